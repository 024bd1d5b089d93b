// TDVP linear solve and time integration on the device (FP64, one CTA):
// SolveForParametersDot (TDVMC.cpp:1713-1828) with the system of
// BuildSystemOfEquationsForParametersIncludePhi (TDVMC.cpp:1506-1537), the
// diagonal preconditioning (1684-1701), the regularisation (1703-1711), the
// Cholesky factorisation and solves (1560-1622) or a pivoted dense solve with
// the mean of the solution removed (type 1, 1763-1827), CalculatePhiDot
// (1658-1682), and the Euler / RK4 / predictor-corrector parameter updates
// (1834-1858, 1969-2035, 1912-1967)
// with NormalizeWavefunction (2525-2529).
//
// Stage bookkeeping lives in DynState so the same captured graph serves all
// four RK4 stages: the kernel reads `stage`, writes the stage derivative and
// the parameters of the next sampling pass, and advances `stage` and the
// Philox `pass` counter.
#pragma once

#include "common.cuh"

namespace tdvmc {

struct SolveArgs {
	int p;
	int imag;        // IMAGINARY_TIME
	int precond;     // USE_PRECONDITIONING
	int solver;      // LINEAR_EQUATION_SOLVER_TYPE (0 Cholesky, 1 pivoted dense)
	int mode;        // 0: right-hand side only, 1: RK4 stage, 2: Euler step, 3: predictor-corrector stage
	int normalize;   // USE_NORMALIZE_WF
	int ldS, ldC;    // leading dimensions of S and of the covariance rows
	int adj_force;   // imaginary time: add half the walker mean of dE_loc/d uR to the force
	int dE_col;      // column of Re dE_loc/d uR_0 in means1 (pairs Re, Im per parameter)
	double dt;
};

// Corrector passes of the predictor-corrector on stored samples (PCsteps in
// CalculateNextParametersPCReuseSamples, TDVMC.cpp:1912-1967): stage 0 is the
// Euler predictor u + u'(u) dt, stage c = 1..kPcCorrectors sets
// u + (u'(u) + u'(trial)) dt / 2 and the last one ends the step.
constexpr int kPcCorrectors = 6;

constexpr int kStatusNotPD = 1;
constexpr int kStatusNonFinite = 2;

// The solve and stage update of one system by one CTA (dynamic shared memory:
// solve_smem_bytes(p)).
template <typename T>
__device__ __forceinline__ void solve_stage(SolveArgs a, DynState* __restrict__ dyn, const double* __restrict__ means1,
                                            const double* __restrict__ S, const double* __restrict__ cov,
                                            const T* __restrict__ lnpsi_w, double* __restrict__ base,
                                            double* __restrict__ stage_params, double* __restrict__ kdot,
                                            double* __restrict__ rhs_out, double* __restrict__ means_step0,
                                            int n_means) {
	extern __shared__ double sm[];
	const int P = a.p;
	const int np = 2 * P + 2;
	double* M = sm;                 // P*(P+2): matrix with two right-hand-side columns
	double* sc = M + P * (P + 2);   // P scales
	double* od = sc + P;            // P original diagonal
	double* sol = od + P;           // 2P solutions (R then I)
	double* tmp = sol + 2 * P;      // 2P
	__shared__ int bad;
	__shared__ int stage_s;
	const int tid = threadIdx.x;
	const int ld = P + 2;
	if (tid == 0) {
		bad = 0;
		stage_s = (a.mode == 1 || a.mode == 3) ? (int)dyn->stage : 0;
	}
	const double* Om = means1;       // <O_k>
	const double ER = means1[P];
	const double EI = means1[P + 1];
	for (int e = tid; e < P * P; e += blockDim.x) {
		const int i = e / P, j = e % P;
		M[i * ld + j] = S[(size_t)i * a.ldS + j];
	}
	for (int i = tid; i < P; i += blockDim.x) {
		const double cR = cov[(size_t)i * a.ldC + 0];  // cov(O_i, E^R)
		const double cI = cov[(size_t)i * a.ldC + 1];  // cov(O_i, E^I)
		double fr, fi;
		if (a.imag == 0) {
			fr = cI;   // <O E^I> - <E^I><O>
			fi = -cR;  // -<O E^R> + <E^R><O>
		} else {
			fr = -cR;
			fi = -(cI + Om[i] * EI);  // -<O E^I>, not centred in the reference
			// adjoint-driven ground-state preparation: -1/2 d<E>/d uR_k with
			// d<E>/d uR_k = 2 cov(O_k, E^R) + <dE_loc/d uR_k>
			if (a.adj_force) fr -= 0.5 * means1[a.dE_col + 2 * i];
		}
		M[i * ld + P] = fr;
		M[i * ld + P + 1] = fi;
	}
	__syncthreads();
	if (a.precond) {
		for (int i = tid; i < P; i += blockDim.x) sc[i] = sqrt(M[i * ld + i]);
		__syncthreads();
		for (int e = tid; e < P * (P + 2); e += blockDim.x) {
			const int i = e / ld, j = e % ld;
			M[e] = (j < P) ? M[e] / (sc[i] * sc[j]) : M[e] / sc[i];
		}
		__syncthreads();
	}
	const double eps = (a.solver == 0) ? 1e-3 : (a.precond ? 2e-3 : 0.0);
	for (int i = tid; i < P; i += blockDim.x) {
		M[i * ld + i] += eps;
		od[i] = M[i * ld + i];
	}
	__syncthreads();

	if (a.solver == 0) {
		// right-looking Cholesky of the lower triangle; a non-positive pivot keeps
		// the original diagonal entry and flags the step, as the reference does
		for (int j = 0; j < P; j++) {
			if (tid == 0) {
				const double d = M[j * ld + j];
				if (d > 0) M[j * ld + j] = sqrt(d);
				else {
					M[j * ld + j] = od[j];
					bad = 1;
				}
			}
			__syncthreads();
			for (int i = j + 1 + tid; i < P; i += blockDim.x) M[i * ld + j] /= M[j * ld + j];
			__syncthreads();
			const int m = P - j - 1;
			for (int e = tid; e < m * m; e += blockDim.x) {
				const int i = j + 1 + e / m, k = j + 1 + e % m;
				if (k <= i) M[i * ld + k] -= M[i * ld + j] * M[k * ld + j];
			}
			__syncthreads();
		}
		// forward / backward substitution: warp 0 -> real rhs, warp 1 -> imaginary rhs
		const int wid = tid >> 5, lane = tid & 31;
		if (wid < 2) {
			const int col = P + wid;
			for (int i = 0; i < P; i++) {
				double s = 0.0;
				for (int j = lane; j < i; j += 32) s += M[i * ld + j] * tmp[wid * P + j];
				for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
				if (lane == 0) tmp[wid * P + i] = 1.0 / M[i * ld + i] * (M[i * ld + col] - s);
				__syncwarp();
			}
			for (int i = P - 1; i >= 0; i--) {
				double s = 0.0;
				for (int j = i + 1 + lane; j < P; j += 32) s += M[j * ld + i] * sol[wid * P + j];
				for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
				if (lane == 0) sol[wid * P + i] = 1.0 / M[i * ld + i] * (tmp[wid * P + i] - s);
				__syncwarp();
			}
		}
		__syncthreads();
	} else {
		// Gaussian elimination with partial pivoting on [M | rhs_R rhs_I]
		__shared__ int piv;
		for (int c = 0; c < P; c++) {
			if (tid == 0) {
				int pv = c;
				for (int r = c + 1; r < P; r++)
					if (fabs(M[r * ld + c]) > fabs(M[pv * ld + c])) pv = r;
				piv = pv;
			}
			__syncthreads();
			if (piv != c)
				for (int j = tid; j < ld; j += blockDim.x) {
					const double t = M[c * ld + j];
					M[c * ld + j] = M[piv * ld + j];
					M[piv * ld + j] = t;
				}
			__syncthreads();
			const int m = P - c - 1;
			for (int e = tid; e < m * (ld - c); e += blockDim.x) {
				const int r = c + 1 + e / (ld - c), j = c + e % (ld - c);
				if (j == c) continue;
				M[r * ld + j] -= M[r * ld + c] / M[c * ld + c] * M[c * ld + j];
			}
			__syncthreads();
			for (int r = c + 1 + tid; r < P; r += blockDim.x) M[r * ld + c] = 0.0;
			__syncthreads();
		}
		const int wid = tid >> 5, lane = tid & 31;
		if (wid < 2) {
			const int col = P + wid;
			for (int i = P - 1; i >= 0; i--) {
				double s = 0.0;
				for (int j = i + 1 + lane; j < P; j += 32) s += M[i * ld + j] * sol[wid * P + j];
				for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
				if (lane == 0) sol[wid * P + i] = (M[i * ld + col] - s) / M[i * ld + i];
				__syncwarp();
			}
			// remove the mean of the solution vector (TDVMC.cpp:1802-1809)
			double s = 0.0;
			for (int j = lane; j < P; j += 32) s += sol[wid * P + j];
			for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
			const double mean = s / P;
			for (int j = lane; j < P; j += 32) sol[wid * P + j] -= mean;
		}
		__syncthreads();
	}

	if (tid == 0) {
		// CalculatePhiDot before the preconditioning scale is undone (as the reference)
		double pr = 0.0, pi = 0.0;
		for (int i = 0; i < P; i++) {
			pr -= Om[i] * sol[i];
			pi -= Om[i] * sol[P + i];
		}
		if (a.imag == 0) pi -= ER;
		else pr -= ER;
		tmp[0] = pr;
		tmp[1] = pi;
	}
	__syncthreads();
	const double phiDotR = tmp[0], phiDotI = tmp[1];
	const int stage = stage_s;
	// slot of this stage's derivative: RK4 one per stage; predictor-corrector: the
	// predictor's in slot 0, the latest corrector's in slot 1
	double* kd = kdot + (size_t)(a.mode == 3 ? (stage == 0 ? 0 : 1) : stage) * np;
	for (int i = tid; i < P; i += blockDim.x) {
		double r = sol[i], im = sol[P + i];
		if (a.precond) {
			r /= sc[i];
			im /= sc[i];
		}
		kd[i] = r;
		kd[P + i] = im;
		if (a.mode == 0) {
			rhs_out[i] = r;
			rhs_out[P + i] = im;
		}
	}
	if (tid == 0) {
		kd[2 * P] = phiDotR;
		kd[2 * P + 1] = phiDotI;
		if (a.mode == 0) {
			rhs_out[2 * P] = phiDotR;
			rhs_out[2 * P + 1] = phiDotI;
		}
	}
	if ((a.mode == 1 || a.mode == 3) && stage == 0)
		for (int i = tid; i < n_means; i += blockDim.x) means_step0[i] = means1[i];
	__syncthreads();

	if (a.mode == 0) {
		if (tid == 0) {
			int st = bad ? kStatusNotPD : 0;
			for (int i = 0; i < np; i++)
				if (!isfinite(rhs_out[i])) st |= kStatusNonFinite;
			dyn->status |= st;
		}
		return;
	}
	const bool last = a.mode == 2 || (a.mode == 1 && stage == 3) || (a.mode == 3 && stage == kPcCorrectors);
	if (last) {
		// final update of the step
		for (int i = tid; i < np; i += blockDim.x) {
			double inc;
			if (a.mode == 2) inc = kdot[i];
			else if (a.mode == 3) inc = (kdot[i] + kdot[np + i]) / 2.0;
			else inc = (kdot[i] + 2.0 * kdot[np + i] + 2.0 * kdot[2 * np + i] + kdot[3 * np + i]) / 6.0;
			base[i] = base[i] + inc * a.dt;
		}
		__syncthreads();
		if (tid == 0 && a.normalize) base[2 * P] = -(double)lnpsi_w[0];
		__syncthreads();
		for (int i = tid; i < np; i += blockDim.x) stage_params[i] = base[i];
	} else if (a.mode == 3) {
		// the predictor, or the next corrector's trial parameters
		for (int i = tid; i < np; i += blockDim.x)
			stage_params[i] = stage == 0 ? base[i] + kdot[i] * a.dt : base[i] + (kdot[i] + kdot[np + i]) * (a.dt / 2.0);
	} else {
		const double cdt = (stage < 2) ? a.dt / 2.0 : a.dt;
		for (int i = tid; i < np; i += blockDim.x) stage_params[i] = base[i] + kd[i] * cdt;
	}
	__syncthreads();
	if (tid == 0) {
		int st = 0;
		if (bad) st |= kStatusNotPD;
		for (int i = 0; i < np; i++)
			if (!isfinite(stage_params[i])) st |= kStatusNonFinite;
		dyn->status |= st;
		dyn->stage = ((a.mode == 1 && stage < 3) || (a.mode == 3 && stage < kPcCorrectors)) ? (uint32_t)(stage + 1) : 0u;
		dyn->pass += 1u;
	}
}

template <typename T>
__global__ void __launch_bounds__(256) k_solve(SolveArgs a, DynState* __restrict__ dyn, const double* __restrict__ means1,
                                               const double* __restrict__ S, const double* __restrict__ cov,
                                               const T* __restrict__ lnpsi_w, double* __restrict__ base,
                                               double* __restrict__ stage_params, double* __restrict__ kdot,
                                               double* __restrict__ rhs_out, double* __restrict__ means_step0,
                                               int n_means) {
	solve_stage<T>(a, dyn, means1, S, cov, lnpsi_w, base, stage_params, kdot, rhs_out, means_step0, n_means);
}

// Independent systems, one CTA each (system b = blockIdx.x): its state, means
// (n_means per system), S (p x p), covariances (p x 2), walkers (nws per
// system, the first one normalises), parameter vectors (2p + 2 per system; the
// RK slopes 4 x (2p + 2)).
template <typename T>
__global__ void __launch_bounds__(256) k_solve_systems(SolveArgs a, DynState* __restrict__ dyn,
                                                       const double* __restrict__ means1, const double* __restrict__ S,
                                                       const double* __restrict__ cov, const T* __restrict__ lnpsi_w,
                                                       int64_t nws, double* __restrict__ base,
                                                       double* __restrict__ stage_params, double* __restrict__ kdot,
                                                       double* __restrict__ rhs_out, double* __restrict__ means_step0,
                                                       int n_means) {
	const size_t b = blockIdx.x;
	const size_t np = 2 * (size_t)a.p + 2;
	solve_stage<T>(a, dyn + b, means1 + b * n_means, S + b * a.p * a.p, cov + b * a.p * 2, lnpsi_w + b * nws,
	               base + b * np, stage_params + b * np, kdot + b * 4 * np, rhs_out + b * np,
	               means_step0 + b * n_means, n_means);
}

__host__ __device__ inline size_t solve_smem_bytes(int p) { return ((size_t)p * (p + 2) + 6 * (size_t)p + 8) * sizeof(double); }

// Stage coefficient tables from the current stage parameters: per-spline
// complex weights w_s = sum_k alpha_k fold[k][s], then per knot interval j the
// cubic sum_q w_{j+3-q} loc[j][q][.]: the real cubic for the sampler, the
// first and second r-derivatives of the complex cubic for the evaluation,
// and the outer-pair value uR[p-1].
template <typename T>
__global__ void __launch_bounds__(128) k_prep(int p, int ns, int nbin, int ncoef, int uniform, double hinv,
                                              const T* __restrict__ hv, const double* __restrict__ params,
                                              const double* __restrict__ fold, const double* __restrict__ loc,
                                              T* __restrict__ coefU, T* __restrict__ coefC, T* __restrict__ uout) {
	__shared__ double wR[kMaxSplines], wI[kMaxSplines];
	for (int s = threadIdx.x; s < ns; s += blockDim.x) {
		double r = 0.0, im = 0.0;
		for (int k = 0; k < p; k++) {
			const double f = fold[(size_t)k * ns + s];
			r += params[k] * f;
			im += params[p + k] * f;
		}
		wR[s] = r;
		wI[s] = im;
	}
	__syncthreads();
	for (int j = threadIdx.x; j < nbin; j += blockDim.x) {
		double cr[4] = {0, 0, 0, 0}, ci[4] = {0, 0, 0, 0};
		for (int q = 0; q < 4; q++) {
			const int s = j + 3 - q;
			const double* l = loc + ((size_t)j * 4 + q) * 4;
			for (int c = 0; c < 4; c++) {
				cr[c] += wR[s] * l[c];
				ci[c] += wI[s] * l[c];
			}
		}
		// evaluation table: du/dr = a0 + t (a1 + t a2), d2u/dr2 = b0 + t b1 with
		// the interval's 1/h folded in; per interval three 4-vectors
		// {a0R a1R a2R b0R} {a0I a1I a2I b0I} {b1R b1I 0 0}
		// 1/h as the kernels of type T see it (with the pieces in their coordinate)
		const double hj = uniform ? (double)(T)hinv : (double)hv[j];
		T* e = coefC + (size_t)j * 12;
		e[0] = (T)(cr[1] * hj);
		e[1] = (T)(2.0 * cr[2] * hj);
		e[2] = (T)(3.0 * cr[3] * hj);
		e[3] = (T)(2.0 * cr[2] * hj * hj);
		e[4] = (T)(ci[1] * hj);
		e[5] = (T)(2.0 * ci[2] * hj);
		e[6] = (T)(3.0 * ci[3] * hj);
		e[7] = (T)(2.0 * ci[2] * hj * hj);
		e[8] = (T)(6.0 * cr[3] * hj * hj);
		e[9] = (T)(6.0 * ci[3] * hj * hj);
		e[10] = e[11] = (T)0;
		// sampler table: the real cubic in tau = t - 1/2 (Taylor shift by 1/2)
		coefU[j * 4 + 0] = (T)(cr[0] + 0.5 * cr[1] + 0.25 * cr[2] + 0.125 * cr[3]);
		coefU[j * 4 + 1] = (T)(cr[1] + cr[2] + 0.75 * cr[3]);
		coefU[j * 4 + 2] = (T)(cr[2] + 1.5 * cr[3]);
		coefU[j * 4 + 3] = (T)cr[3];
	}
	if (threadIdx.x == 0) *uout = (T)params[p - 1];
	// entries nbin.. of the sampler table: the constant outer-pair value
	for (int j = nbin + threadIdx.x; j < ncoef; j += blockDim.x) {
		coefU[j * 4 + 0] = (T)params[p - 1];
		coefU[j * 4 + 1] = coefU[j * 4 + 2] = coefU[j * 4 + 3] = (T)0;
	}
}

}  // namespace tdvmc
