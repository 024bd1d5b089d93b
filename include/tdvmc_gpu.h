/*
 * tdvmc_gpu.h -- C ABI of the GB300 (sm_103a) TDVP hot path.
 *
 * Drop-in for the batched form of the reference's physics plugin and TDVP
 * driver step (mathiasgartner/TDVMC):
 *   - PhysicalSystems::IPhysicalSystem (src/PhysicalSystems/IPhysicalSystem.h:16-123)
 *     as implemented by PhysicalSystems::BosonsBulk
 *     (src/PhysicalSystems/BosonsBulk.cpp), evaluated for all walkers at once;
 *   - the sampling loop DoMetropolisStep / UpdateExpectationValues
 *     (src/TDVMC.cpp:858-924, 1038-1150);
 *   - the rank reduction ParallelUpdateExpectationValues (src/TDVMC.cpp:1152-1220,
 *     src/MPIMethods.h:191-206), here one on-device reduction;
 *   - SolveForParametersDot and the RK4 integrator (src/TDVMC.cpp:1506-1828,
 *     1969-2035).
 *
 * Conventions: every entry point returns an int status (TDVMC_OK = 0, >0 an
 * error code, see tdvmc_status_string); no C++ exception crosses the ABI.
 * Array arguments are HOST pointers with the layouts documented per call;
 * they are copied to/from device memory on the context's CUDA stream and the
 * call returns after the copy-out completes.  A context is bound to the
 * current CUDA device at creation, owns one stream, and is not thread-safe.
 *
 * Walker layout: walker-major structure of arrays, x[w][d][i] for walker w,
 * Cartesian component d < dim and particle i < n (doubles on the host; the
 * device keeps them in the context precision).
 */
#ifndef TDVMC_GPU_H
#define TDVMC_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TDVMC_OK 0
#define TDVMC_ERR_ARG 1        /* invalid argument or size */
#define TDVMC_ERR_CUDA 2       /* a CUDA runtime call failed */
#define TDVMC_ERR_NOMEM 3      /* device allocation failed */
#define TDVMC_ERR_STATE 4      /* call order (e.g. no walkers set) */
#define TDVMC_ERR_NOT_PD 5     /* Cholesky met a non-positive pivot (reference: doNotAcceptStep) */
#define TDVMC_ERR_NONFINITE 6  /* a non-finite parameter or energy was produced */

/* arithmetic of the walker / pair kernels */
#define TDVMC_PREC_FP64 0  /* plain FP64 everywhere */
#define TDVMC_PREC_MIXED 1 /* FP32 pairs and walkers, 3xTF32 tensor-core S, FP64 centring/solve/RK4 */

/* pair potentials; parameters [a, b, t_quench, a', b'] as BosonsBulk.cpp:237-242 */
#define TDVMC_POT_NONE 0
#define TDVMC_POT_SQUARE 1 /* b if r < a           (BosonsBulk.cpp:268-271) */
#define TDVMC_POT_GAUSS 2  /* b exp(-(r/a)^2 / 2)  (BosonsBulk.cpp:263-265)  */
#define TDVMC_POT_LJ 3     /* 4 b ((a/r)^12 - (a/r)^6) (Potentials/LJ.cpp:16-22) */

/* physical systems: the reference's SYSTEM_TYPE (src/TDVMC.cpp:2843-2850, 2953-2960) */
#define TDVMC_SYS_BOSONS_BULK 0 /* PhysicalSystems::BosonsBulk */
/* PhysicalSystems::NUBosonsBulkPB: a pair at r >= r_max enters every sum at the
 * mirrored distance r' = 2 r_max - r and counts iff r' < r_max; gradient terms
 * d / r' with the sign of d (NUBosonsBulkPB.cpp:333-336, 381-392); Laplacian
 * (D-1)/r' (398); square-well potential b [r' < a] (347-350); boundary fold
 * O_k = S_{k+1}, O_1 += S_0, O_{p-1} += S_{p+1} (219-228).  Requires the knots
 * (n_user_knots = p: the reference reads them before it builds any default),
 * pot_kind TDVMC_POT_SQUARE, and 2 r_max >= sqrt(dim) L / 2 so that every
 * mirrored distance is non-negative (below that the reference indexes its
 * spline tables out of range). */
#define TDVMC_SYS_NU_BOSONS_BULK_PB 1
/* NUBosonsBulkPB with the exact derivatives of the mirrored pair term
 * u(2 r_max - r): at a pair beyond r_max the gradient term is -u'(r') d / r and
 * the Laplacian's -(D-1)/r u'(r') (d r'/d r = -1, the sign flip the reference
 * has commented out at NUBosonsBulkPB.cpp:387); ln psi, O_k, the moves and the
 * potential as TDVMC_SYS_NU_BOSONS_BULK_PB. */
#define TDVMC_SYS_NU_BOSONS_BULK_PB_EXACT 2

typedef struct tdvmc_ctx tdvmc_ctx;

/* System description: the reference's globals N, DIM, N_PARAM, LBOX
 * (src/TDVMC.cpp:84-89), SYSTEM_PARAMS, NURBS_GRID (TDVMC.cpp:128-131),
 * SYSTEM_TYPE and the compile-time HBAR2_2M (src/Constants.h:12), plus the
 * walker count.  Zero-initialise it (`tdvmc_system_desc d = {};`): a field
 * left 0 takes its default (system_type 0 is BosonsBulk). */
typedef struct tdvmc_system_desc {
	int32_t dim;               /* 1, 2 or 3 */
	int32_t n;                 /* particles per walker, 2..1024 */
	int32_t p;                 /* variational parameters (N_PARAM), 4..128 */
	int32_t n_user_knots;      /* 0: uniform knots on [0, L/2] (BosonsBulk.cpp:61-67) */
	const double* user_knots;  /* n_user_knots values (SetNodes, BosonsBulk.cpp:35-44); must equal p */
	double box_length;         /* LBOX */
	int32_t pot_kind;          /* TDVMC_POT_* */
	int32_t n_pot;             /* number of entries used in pot[] (2 or 5) */
	double pot[5];
	double hbar2_2m;           /* HBAR2_2M; 1.0 in the reference */
	int32_t precision;         /* TDVMC_PREC_* */
	int32_t system_type;       /* TDVMC_SYS_*; 0 (zero-initialised) is BosonsBulk */
	int64_t n_walkers;         /* independent Markov chains, >= 1 */
} tdvmc_system_desc;

/* Walker-mean statistics of the last evaluation, FP64.  The moments are the
 * reference's accumulators (TDVMC.cpp:147-153) after ReduceToAverage, with S
 * and the force already centred (S_kl = <O_k O_l> - <O_k><O_l>). */
typedef struct tdvmc_stats {
	int64_t n_walkers;
	double energy_re, energy_im;   /* <E^R>, <E^I> */
	double other[9];               /* otherExpectationValues (BosonsBulk.cpp:449-457) */
	double accept_rate;            /* accepted / proposed moves of the last sampling pass */
	int32_t status;                /* TDVMC_OK or TDVMC_ERR_NOT_PD / NONFINITE of the last solve */
	int32_t reserved;
} tdvmc_stats;

/* Options of one TDVP step. */
typedef struct tdvmc_step_opts {
	double dt;                 /* TIMESTEP */
	int32_t imaginary_time;    /* IMAGINARY_TIME: 0 real, 1 imaginary */
	int32_t ode_solver;        /* ODE_SOLVER_TYPE: 0 Euler, 2 RK4, 3 RK4 on stored samples,
	                              5 predictor-corrector on stored samples (Euler predictor,
	                              6 trapezoidal corrector passes, CalculateNextParametersPCReuseSamples) */
	int32_t lin_solver;        /* LINEAR_EQUATION_SOLVER_TYPE: 0 Cholesky (+1e-3 I) */
	int32_t precondition;      /* USE_PRECONDITIONING */
	int32_t normalize_wf;      /* USE_NORMALIZE_WF: phiR <- -ln psi of walker 0 */
	int32_t moves_per_stage;   /* single-particle moves per walker per sampling pass (MC_NTHERMSTEPS) */
	double mc_step;            /* MC_STEP: Gaussian displacement width */
	uint64_t seed;             /* Philox key */
	int32_t use_adjoint;       /* 1: also compute <dE_loc/d alpha> each stage; 2: in imaginary time
	                              also drive the force with it, F_k = -(cov(O_k, E^R) + <dE_loc/d uR_k>/2),
	                              i.e. -1/2 d<E>/d uR_k (no reference counterpart) */
	int32_t update_every;      /* ode_solver 3, 5: UPDATE_SAMPLES_EVERY_NTH_STEP; 0 samples every walker each step,
	                              k > 0 refreshes a window of walkers every k-th step */
	double update_percent;     /* ode_solver 3, 5: UPDATE_SAMPLES_PERCENT, size of the refresh window in % of walkers */
} tdvmc_step_opts;

const char* tdvmc_status_string(int status);

/* Create / destroy.  Replaces IPhysicalSystem construction + InitSystem
 * (BosonsBulk.cpp:8-156) for n_walkers walkers.  Fails with TDVMC_ERR_ARG
 * on the parameter-count mismatch that makes the reference exit
 * (BosonsBulk.cpp:85-91). */
int tdvmc_create(const tdvmc_system_desc* desc, tdvmc_ctx** out);
int tdvmc_destroy(tdvmc_ctx* ctx);
/* the context's CUDA stream (cudaStream_t), for callers that time or order work */
int tdvmc_get_stream(tdvmc_ctx* ctx, void** stream);

/* IPhysicalSystem::SetTime (IPhysicalSystem.h:70): selects the quench branch
 * of the pair potential (BosonsBulk.cpp:239-242). */
int tdvmc_set_time(tdvmc_ctx* ctx, double time);

/* Parameters uR[p], uI[p], phiR, phiI (BroadcastNewParameters, TDVMC.cpp:506-512). */
int tdvmc_set_params(tdvmc_ctx* ctx, const double* uR, const double* uI, double phiR, double phiI);
int tdvmc_get_params(tdvmc_ctx* ctx, double* uR, double* uI, double* phiR, double* phiI);

/* Walker coordinates, layout x[w][d][i] (nw = n_walkers). */
int tdvmc_set_walkers(tdvmc_ctx* ctx, const double* x, int64_t nw);
int tdvmc_get_walkers(tdvmc_ctx* ctx, double* x, int64_t nw);

/* `moves` single-particle Metropolis moves per walker (DoMetropolisStep,
 * TDVMC.cpp:858-916) with the current parameters.  Random numbers: Philox
 * with key `seed` and counter {move, walker, pass, call}.  *accepted (may be
 * NULL) receives the total number of accepted moves. */
int tdvmc_sample(tdvmc_ctx* ctx, int32_t moves, double mc_step, uint64_t seed, uint32_t pass, int64_t* accepted);

/* Forward evaluation at the current walkers (CalculateWavefunction +
 * CalculateExpectationValues, BosonsBulk.cpp:179-545).  Outputs (any may be
 * NULL): lnpsi[nw]; O[nw*p] walker-major; eloc[nw*2] = (E^R, E^I);
 * other7[nw*7] = {kineticR, V_int, sumR1, sumI1, sumR2, sumI2, sumR1I1}.
 * The first evaluation of a context allocates its particle-gradient scratch
 * (nw x 6 x n values; TDVMC_ERR_NOMEM if it does not fit), which the forward
 * and adjoint sweeps share. */
int tdvmc_eval_local(tdvmc_ctx* ctx, double* lnpsi, double* O, double* eloc, double* other7);

/* Backward: the same forward pass plus one reverse sweep over the pairs,
 * giving dE[nw*p*2] = (Re, Im) of dE_loc/d uR_k (holomorphic: d/d uI_k is
 * i times it).  Minimum-image distances are recomputed, no pair table is
 * stored.  No counterpart exists in the reference (its force is the SR
 * covariance only, TDVMC.cpp:1527-1528). */
int tdvmc_eval_local_adjoint(tdvmc_ctx* ctx, double* dE);

/* Correlated sampling.  tdvmc_store_samples keeps, for every walker at its
 * current position, the parameter-independent data of the local quantities
 * (InitCorrelatedSamplingData + FillCorrelatedSamplingData,
 * BosonsBulk.cpp:667-681; CSDataBulkSplines.h:9-16): per spline and particle
 * sum_i B'(r) rhat, the summed B'' + (D-1)/r B', O_k, V_int and the outer-pair
 * count.  nw * (p+2) * 3 * n32 values of the working precision, n32 = n
 * rounded up to a multiple of 32 (8.9 GB in FP32 at nw = 65,536, n = 343,
 * p = 30); the store is allocated on first use (TDVMC_ERR_NOMEM if it does
 * not fit).
 * Moving the walkers (tdvmc_set_walkers, tdvmc_sample, a resampling step)
 * invalidates it. */
int tdvmc_store_samples(tdvmc_ctx* ctx);

/* Local quantities of the stored samples at the current parameters, without
 * resampling (CalculateWavefunction + CalculateExpectationValues for an
 * ICorrelatedSamplingData, BosonsBulk.cpp:468-472, 547-551).  Same outputs
 * as tdvmc_eval_local, plus dE as tdvmc_eval_local_adjoint when dE is not
 * NULL.  ln psi uses the sample's own outer-pair count (the reference uses
 * that of the configuration it evaluated last).  TDVMC_ERR_STATE without a
 * valid store. */
int tdvmc_eval_stored(tdvmc_ctx* ctx, double* lnpsi, double* O, double* eloc, double* other7, double* dE);

/* Pair distribution and static structure factor of the current walkers,
 * averaged over walkers (BosonsBulk::CalculateAdditionalSystemProperties,
 * BosonsBulk.cpp:474-520; each walker is one sample of the running mean of
 * CalculateAdditionalSystemProperties, TDVMC.cpp:1332-1388).
 * g(r): the grid [0, r_max) with spacing r_max / gr_bins (GR_BIN_COUNT,
 * BosonsBulk.cpp:145); gr[] receives *gr_count (<= gr_bins) values: pairs
 * i < j with r < r_max, each adding D/(N-1) / (volume of its shell)
 * (NUBosonsBulkPB: 1 / (volume of its shell), NUBosonsBulkPB.cpp:602-612).
 * S(k): kvec[nvec*dim] are the k vectors already scaled by 2 pi / L (the
 * integer vectors of kVectors{D}D.json), shell s owns rows
 * shell_off[s] .. shell_off[s+1]-1 (shell_off[0] = 0, nvec <= 4096);
 * sk[s] = |sum over the shell's vectors and the particles of exp(i k.r)|^2 /
 * (N * vectors in the shell).  nshell = 0 skips S(k). */
int tdvmc_observables(tdvmc_ctx* ctx, int32_t gr_bins, int32_t nshell, const int32_t* shell_off, const double* kvec,
                      double* gr, int32_t* gr_count, double* sk);

/* Walker-mean reduction of the last evaluation (ParallelUpdateExpectationValues,
 * TDVMC.cpp:1152-1220).  Optional outputs: O_mean[p], S[p*p] (centred),
 * cov_OER[p], cov_OEI[p], dE_mean[2p] (zeros unless the last evaluation was
 * the adjoint one). */
int tdvmc_reduce_stats(tdvmc_ctx* ctx, tdvmc_stats* stats, double* O_mean, double* S, double* cov_OER,
                       double* cov_OEI, double* dE_mean);

/* SolveForParametersDot (TDVMC.cpp:1713-1828) on the last reduction.
 * Returns TDVMC_ERR_NOT_PD (with the outputs filled as the reference would)
 * when the Cholesky met a non-positive pivot. */
int tdvmc_tdvp_rhs(tdvmc_ctx* ctx, int32_t imaginary_time, int32_t precondition, int32_t lin_solver,
                   double* uDotR, double* uDotI, double* phiDotR, double* phiDotI);

/* One TDVP time step (CalculateNextParameters with ODE_SOLVER_TYPE 0 or 2,
 * TDVMC.cpp:1834-1858, 1969-2035, including the stage-1 sampling of the main
 * loop, TDVMC.cpp:3656): each stage is one CUDA-graph launch of
 * sample -> evaluate (+adjoint) -> reduce -> solve.  Parameters are updated
 * on the device; `stats` (may be NULL) receives the statistics of the first
 * stage, which the reference records per step (TDVMC.cpp:3748-3755).  The
 * Philox pass counter advances by one per stage. */
int tdvmc_step(tdvmc_ctx* ctx, const tdvmc_step_opts* opts, tdvmc_stats* stats);

/* Walker means <O_k> (p values) and the FP64 means of the first stage of the
 * last step (the localOperators the reference records per step,
 * TDVMC.cpp:3750). */
int tdvmc_get_step_operators(tdvmc_ctx* ctx, double* O_mean);

/* `nsteps` steps back to back without host synchronisation (benchmarking
 * and long runs); statistics of the last step's first stage in *stats. */
int tdvmc_run_steps(tdvmc_ctx* ctx, const tdvmc_step_opts* opts, int32_t nsteps, tdvmc_stats* stats);

/* Run `nsteps` steps as tdvmc_run_steps and return the device time between
 * two CUDA events recorded on the context stream around them (*ms).  For
 * benchmarking; no reference counterpart (the reference times whole steps
 * on the host, TDVMC.cpp:3400-3423). */
int tdvmc_time_steps(tdvmc_ctx* ctx, const tdvmc_step_opts* opts, int32_t nsteps, float* ms);

/* Run ONE stage of a step eagerly (no graph) with a CUDA event pair around
 * every kernel; ms[i] receives the duration of kernel i and names[i] (may be
 * NULL) a static name.  *count receives the number of kernels (<= 16).
 * The stage moves the walkers and the Philox pass counter like a graph launch
 * would; the parameters and the stage index are then put back to the step
 * boundary the call started from (base parameters, stage 0), so that the next
 * step is a whole step. */
int tdvmc_profile_stage(tdvmc_ctx* ctx, const tdvmc_step_opts* opts, float* ms, const char** names, int32_t* count);

/* Choose the group width (lanes per walker) and walkers per block of the
 * sampling and evaluation kernels by timing the candidates on the current
 * walkers.  Results are kept in the context. */
int tdvmc_autotune(tdvmc_ctx* ctx, int32_t moves, double mc_step);
/* Report the chosen tiles: lanes per walker and walkers per block of the
 * sampler and the evaluation kernels (evaluation walkers per block 0: each
 * evaluation kernel takes the count in {1, 2, 4} that keeps the most walkers
 * resident per SM). */
int tdvmc_get_tiles(tdvmc_ctx* ctx, int32_t* sample_lanes, int32_t* sample_walkers_per_block,
                    int32_t* eval_lanes, int32_t* eval_walkers_per_block);

/* Measurement utility: FP32 FMA throughput of the current device in
 * TFLOP/s (dependent-free FMA loop on every SM), the ceiling of the
 * CUDA-core-bound sampling and evaluation kernels.  No reference counterpart. */
int tdvmc_measure_fp32_peak(double* tflops);

/* Walker statistics without any device allocation.
 *
 * For callers that cannot allocate device memory, e.g. a host program that
 * owns all GPU memory through its own pool allocator and forbids cudaMalloc /
 * cudaFree while it runs: they pass device arrays they already own.  Computes
 * from O[nw*p] (walker-major) and eloc[nw*2] (E^R, E^I) the same FP64 results
 * as tdvmc_reduce_stats: O_mean[p], E_mean[2], the centred S[p*p] and
 * cov_OER[p], cov_OEI[p].  All pointers are device pointers; the work is
 * queued on `stream` (a cudaStream_t, NULL for the default stream) and the
 * call returns without waiting for it.
 *
 * Limit: p <= 32.  Larger p returns TDVMC_ERR_ARG.  The partial sums live in
 * one fixed file-scope device array of about 0.6 MB that every device which
 * loads this library keeps until the process exits; the call itself
 * allocates nothing.  The first call on a device looks up that array's
 * device address with the device current, so make the first call on each
 * device before any stream capture.  All calls share the array: calls whose
 * work overlaps on the GPU (other streams or host threads) race on it.  A CUDA
 * error already pending on the calling thread is left in place and returned
 * as TDVMC_ERR_CUDA without launching anything.
 *
 * No counterpart in the reference (its averages live in host vectors,
 * TDVMC.cpp:1103-1109). */
int tdvmc_reduce_walkers_noalloc(const double* O, const double* eloc, int64_t nw, int32_t p, double* O_mean,
                                 double* E_mean, double* S, double* cov_OER, double* cov_OEI, void* stream);

/* Number of kernel launches issued by this context since creation. */
int64_t tdvmc_launch_count(tdvmc_ctx* ctx);

/* ------------------------------------------------------------------------
 * Batched trapped drops: many independent 3D systems of uneven particle
 * number, each with its own parameters, walkers, statistics and TDVP solve,
 * every kernel one launch over all drops (persistent blocks taking work items
 * of one drop from a device queue, drops with more particles first).
 *
 * A drop of n bosons (2..32) has open boundaries and
 *   ln psi = sum_k alpha_k O_k + alpha_p sum_i |r_i|^2 + phi,
 * where O_k (k < p) are the BC-folded pair-spline sums of BosonsBulk on
 * uniform knots over [0, r_max] (with its outer-pair term alpha_{p-1} for
 * pairs beyond r_max, BosonsBulk.cpp:61-87, 179-218, 522-545), evaluated with
 * plain displacements as the open-boundary cluster systems do
 * (BosonCluster.cpp:14 USE_NIC = false), and O_p = sum_i |r_i|^2 is the
 * one-body Gaussian width.  Potential: the harmonic trap
 * omega^2 / (4 hbar2_2m) |r|^2 ((m/2) omega^2 r^2 with hbar = 1) plus the
 * Gaussian pair repulsion v0 exp(-r^2 / (2 sigma^2)) over all pairs.  No
 * reference system has this form; the pair-spline part is the BosonsBulk
 * algorithm (same fold, kinetic sums, adjoint) without the minimum image.
 * With v0 = 0, alpha_k = 0 (k < p) and alpha_p = -omega / (4 hbar2_2m) the
 * wave function is the exact ground state: E_loc = (3/2) omega n for every
 * configuration.
 *
 * Per-drop arrays are drop-major: parameters [S][p+1], walker outputs
 * [S][walkers][...], walkers x[s][w][d][i] concatenated over drops. */
typedef struct tdvmc_drops tdvmc_drops;

typedef struct tdvmc_drops_desc {
	int32_t n_systems;         /* S >= 1 */
	const int32_t* n;          /* particles per drop, S values in 2..32 */
	int32_t p;                 /* pair-spline parameters per drop, 4..32 (uniform knots) */
	const double* rmax;        /* per drop: range of the pair spline */
	double omega;              /* trap frequency */
	double v0, sigma;          /* Gaussian pair repulsion */
	double hbar2_2m;
	int32_t precision;         /* TDVMC_PREC_* */
	int64_t walkers_per_system;
} tdvmc_drops_desc;

int tdvmc_drops_create(const tdvmc_drops_desc* desc, tdvmc_drops** out);
int tdvmc_drops_destroy(tdvmc_drops* ctx);
int tdvmc_drops_get_stream(tdvmc_drops* ctx, void** stream);
/* uR, uI [S][p+1]; phiR, phiI [S] (either may be NULL: zeros).  Starts a new step. */
int tdvmc_drops_set_params(tdvmc_drops* ctx, const double* uR, const double* uI, const double* phiR,
                           const double* phiI);
int tdvmc_drops_get_params(tdvmc_drops* ctx, double* uR, double* uI, double* phiR, double* phiI);
/* x: S * walkers * 3 * n_s values, x[s][w][d][i]. */
int tdvmc_drops_set_walkers(tdvmc_drops* ctx, const double* x);
int tdvmc_drops_get_walkers(tdvmc_drops* ctx, double* x);
/* moves_per_particle * n_s single-particle moves per walker (DoMetropolisStep,
 * TDVMC.cpp:858-916) at the current parameters; Philox key `seed`, counter
 * {move, s * walkers + w, pass, call}; *accepted: total accepted moves. */
int tdvmc_drops_sample(tdvmc_drops* ctx, int32_t moves_per_particle, double mc_step, uint64_t seed, uint32_t pass,
                       int64_t* accepted);
/* Local quantities of every walker (CalculateWavefunction +
 * CalculateExpectationValues for each drop): lnpsi [S][w], O [S][w][p+1],
 * eloc [S][w][2], other7 [S][w][7] (as tdvmc_eval_local; V = trap + pair),
 * and, when dE is not NULL, the adjoint dE [S][w][p+1][2] (dE_loc/d uR_k,
 * no reference counterpart).  Any output may be NULL. */
int tdvmc_drops_eval(tdvmc_drops* ctx, double* lnpsi, double* O, double* eloc, double* other7, double* dE);
/* Per-drop walker means of the last evaluation (ParallelUpdateExpectationValues,
 * TDVMC.cpp:1152-1220, per drop): O_mean [S][p+1], energy [S][2], centred S
 * [S][p+1][p+1], cov_OER / cov_OEI [S][p+1], dE_mean [S][p+1][2] (zeros
 * without the adjoint), accepted_mean [S] (accepted moves per walker of the
 * last sampling pass).  Any output may be NULL. */
int tdvmc_drops_reduce(tdvmc_drops* ctx, double* O_mean, double* energy, double* S, double* cov_OER,
                       double* cov_OEI, double* dE_mean, double* accepted_mean);
/* SolveForParametersDot (TDVMC.cpp:1713-1828) of every drop on its last
 * reduction: uDotR/uDotI [S][p+1], phiDotR/phiDotI [S], status [S]
 * (TDVMC_OK or TDVMC_ERR_NOT_PD / NONFINITE per drop; may be NULL).  Returns
 * the worst status. */
int tdvmc_drops_tdvp_rhs(tdvmc_drops* ctx, int32_t imaginary_time, int32_t precondition, int32_t lin_solver,
                         double* uDotR, double* uDotI, double* phiDotR, double* phiDotI, int32_t* status);
/* `nsteps` TDVP steps of every drop (ODE_SOLVER_TYPE 0 or 2): each stage is one
 * CUDA-graph launch of prep -> sample -> evaluate (+adjoint) -> per-drop reduce
 * -> per-drop solve.  opts->moves_per_stage is the number of moves PER
 * PARTICLE (sweeps) of a sampling pass.  energy [S][2] (may be NULL): the
 * first-stage energies of the last step; status [S] as tdvmc_drops_tdvp_rhs. */
int tdvmc_drops_run_steps(tdvmc_drops* ctx, const tdvmc_step_opts* opts, int32_t nsteps, double* energy,
                          int32_t* status);
/* The same steps timed with CUDA events on the context stream (*ms). */
int tdvmc_drops_time_steps(tdvmc_drops* ctx, const tdvmc_step_opts* opts, int32_t nsteps, float* ms);
/* One stage eagerly with an event after every kernel (as tdvmc_profile_stage). */
int tdvmc_drops_profile_stage(tdvmc_drops* ctx, const tdvmc_step_opts* opts, float* ms, const char** names,
                              int32_t* count);
/* Choose the walkers per block of the sampling and evaluation kernels from
 * {32, 64, 128} by timing them on the current walkers (restored afterwards). */
int tdvmc_drops_autotune(tdvmc_drops* ctx, int32_t moves_per_particle, double mc_step);
int tdvmc_drops_get_tiles(tdvmc_drops* ctx, int32_t* sample_threads, int32_t* eval_threads);
int64_t tdvmc_drops_launch_count(tdvmc_drops* ctx);

#ifdef __cplusplus
}
#endif
#endif
