// Batched trapped drops: many independent 3D systems of uneven particle
// number in one launch per kernel.  Each drop is a pair-spline Jastrow with
// the BosonsBulk spline machinery (uniform knots on [0, r_max], the boundary
// fold, the outer-pair term uR[p-1] for pairs beyond r_max; BosonsBulk.cpp:
// 61-87, 179-218, 220-336, 349-458, 522-545), open boundaries (plain
// displacements, as the cluster systems: BosonCluster.cpp:14 USE_NIC =
// false), plus one one-body parameter alpha_p with ln psi += alpha_p sum_i
// |r_i|^2, a harmonic trap kappa |r|^2 and a Gaussian pair repulsion
// v0 exp(-r^2 / (2 sigma^2)) over all pairs.
//
// Work is split into items (drop, first walker, walker count); the sampling
// and evaluation kernels are persistent: each block takes the next item from
// a device counter, items ordered by decreasing particle number so that the
// expensive drops start first.  One thread owns one walker: with at most 32
// particles a walker's coordinates, gradients and spline sums fit in a
// thread-private column of shared memory ([row][thread], conflict-free), and
// no cross-lane reduction is needed per move.
#pragma once

#include "common.cuh"
#include "k_sample.cuh"

namespace tdvmc {

constexpr int kDropMaxN = 32;
constexpr int kDropMaxP = 32;  // pair-spline parameters per drop

// Per-drop constants (device table).
struct DropSys {
	int n;           // particles
	int nbin;        // knot intervals on [0, r_max] (p - 1)
	double rmax, hinv;
	float hf, hf_lo;          // 1/h split for the FP32 local coordinate
	float rcut_lo, rcut_hi;   // FP32 band around r_max decided again in FP64
	long long pos_off;        // first coordinate of the drop's walker block
};

// Physics and sizes shared by all drops (kernel parameter).
struct DropConst {
	int p;           // pair-spline parameters; the one-body parameter is index p
	int p1;          // p + 1
	int ns;          // splines p + 2
	int np;          // parameters per drop in the FP64 stage vectors: 2 p1 + 2
	int ncoef;       // sampler table entries per drop (nbin + 1 of the largest drop)
	int nbin_max;    // evaluation table intervals per drop
	int64_t nws;     // walkers per drop
	double v0, inv2s2;  // Gaussian repulsion v0 exp(-r^2 inv2s2)
	double kappa;       // trap coefficient
	double hbar2_2m;
};

// Columns of the per-drop walker means (pass 1 of k_drop_reduce).
struct DropCols {
	int p1;
	__host__ __device__ int ER() const { return p1; }
	__host__ __device__ int EI() const { return p1 + 1; }
	__host__ __device__ int other() const { return p1 + 2; }  // 7
	__host__ __device__ int acc() const { return p1 + 9; }
	__host__ __device__ int dE() const { return p1 + 10; }  // 2 p1
	__host__ __device__ int count() const { return 3 * p1 + 10; }
};

// The next work item of a persistent kernel (block-uniform).
__device__ __forceinline__ int next_item(int* counter) {
	__shared__ int item_s;
	__syncthreads();  // every thread is done with the previous item
	if (threadIdx.x == 0) item_s = atomicAdd(counter, 1);
	__syncthreads();
	return item_s;
}

// Stage tables of every drop from the drop's stage parameters (one block per
// drop): the sampler's real cubic per interval in tau = t - 1/2 plus the
// outer-pair constant, and the evaluation's first and second r-derivatives of
// the complex cubic (layouts of k_prep).  loc[q][c]: the four uniform pieces.
template <typename T>
__global__ void __launch_bounds__(128) k_drop_prep(DropConst dc, const DropSys* __restrict__ sys,
                                                   const double* __restrict__ stage, const double* __restrict__ fold,
                                                   const double* __restrict__ loc, T* __restrict__ coefU,
                                                   T* __restrict__ coefC) {
	__shared__ double wR[kDropMaxP + 2], wI[kDropMaxP + 2];
	const int s = blockIdx.x;
	const DropSys sy = sys[s];
	const double* prm = stage + (size_t)s * dc.np;
	const int P = dc.p, ns = dc.ns, p1 = dc.p1;
	for (int k = threadIdx.x; k < ns; k += blockDim.x) {
		double r = 0.0, im = 0.0;
		for (int q = 0; q < P; q++) {
			const double f = fold[(size_t)q * ns + k];
			r += prm[q] * f;
			im += prm[p1 + q] * f;
		}
		wR[k] = r;
		wI[k] = im;
	}
	__syncthreads();
	T* cu = coefU + (size_t)s * dc.ncoef * 4;
	T* cc = coefC + (size_t)s * dc.nbin_max * 12;
	const double hj = sy.hinv;
	for (int j = threadIdx.x; j < dc.ncoef; j += blockDim.x) {
		if (j >= sy.nbin) {
			cu[j * 4 + 0] = (T)prm[P - 1];
			cu[j * 4 + 1] = cu[j * 4 + 2] = cu[j * 4 + 3] = T(0);
			continue;
		}
		double cr[4] = {0, 0, 0, 0}, ci[4] = {0, 0, 0, 0};
		for (int q = 0; q < 4; q++) {
			const int sp = j + 3 - q;
			for (int c = 0; c < 4; c++) {
				cr[c] += wR[sp] * loc[q * 4 + c];
				ci[c] += wI[sp] * loc[q * 4 + c];
			}
		}
		cu[j * 4 + 0] = (T)(cr[0] + 0.5 * cr[1] + 0.25 * cr[2] + 0.125 * cr[3]);
		cu[j * 4 + 1] = (T)(cr[1] + cr[2] + 0.75 * cr[3]);
		cu[j * 4 + 2] = (T)(cr[2] + 1.5 * cr[3]);
		cu[j * 4 + 3] = (T)cr[3];
		T* e = cc + (size_t)j * 12;
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
		e[10] = e[11] = T(0);
	}
}

// Pair function u(r) of the sampler from r^2 (uniform knots; entries nbin..
// of the table hold the outer-pair constant).
template <typename T>
__device__ __forceinline__ T drop_u(const DropSys& sy, T r2, const Q4<T>* __restrict__ coef) {
	const T r = pair_r(r2);
	const T xm = fma(r, (T)sy.hinv, T(-0.5));
	const T R = sizeof(T) == 4 ? (T)kRoundF : (T)kRoundD;
	T y = xm + R;
	y = fmin(y, R + (T)sy.nbin);
	const T jf = y - R;
	const T tau = xm - jf;
	int j;
	if (sizeof(T) == 4) j = __float_as_int((float)y) - __float_as_int(kRoundF);
	else j = (int)(__double_as_longlong((double)y) - __double_as_longlong(kRoundD));
	const Q4<T> c = coef[j];
	return c.x + tau * (c.y + tau * (c.z + tau * c.w));
}

// Metropolis sampling of every walker of every drop: moves_per_particle * n
// single-particle moves per walker (DoMetropolisStep, TDVMC.cpp:858-916) with
// the direct exponent change sum_i u(r_new) - u(r_old) + alpha_p (|x_new|^2 -
// |x_old|^2); Philox counter {move, global walker, pass, call} as the bulk
// sampler.  Shared memory: the item's table coef[ncoef] | positions
// X[3 nmax][blockDim].
template <typename T>
__global__ void __launch_bounds__(128) k_drop_sample(DropConst dc, const DropSys* __restrict__ sys,
                                                     const int4* __restrict__ items, int nitems,
                                                     int* __restrict__ counter, const T* __restrict__ coefU,
                                                     const double* __restrict__ stage, T* __restrict__ pos,
                                                     int moves_per_particle, T step, uint2 key,
                                                     const DynState* __restrict__ dyn, int nmax,
                                                     int* __restrict__ acc_out) {
	extern __shared__ __align__(32) unsigned char smem_raw[];
	Q4<T>* coef = reinterpret_cast<Q4<T>*>(smem_raw);
	T* X = reinterpret_cast<T*>(coef + dc.ncoef);
	const int tid = threadIdx.x, B = blockDim.x;
	const uint32_t pass = dyn[0].pass;
	for (;;) {
		const int it = next_item(counter);
		if (it >= nitems) break;
		const int4 wi = items[it];
		const int s = wi.x;
		const DropSys sy = sys[s];
		const int n = sy.n;
		for (int i = tid; i < dc.ncoef; i += B) {
			const T* c = coefU + ((size_t)s * dc.ncoef + i) * 4;
			coef[i] = Q4<T>{c[0], c[1], c[2], c[3]};
		}
		const T aP = (T)stage[(size_t)s * dc.np + dc.p];
		__syncthreads();
		if (tid < wi.z) {
			const int64_t w = wi.y + tid;
			const int64_t g = (int64_t)s * dc.nws + w;
			T* pw = pos + sy.pos_off + (size_t)w * 3 * n;
			for (int e = 0; e < 3 * n; e++) X[(size_t)e * B + tid] = pw[e];  // row d*n + i
			const int moves = moves_per_particle * n;
			int nacc = 0;
			for (int m = 0; m < moves; m++) {
				const MoveRand<T> mr = move_rand<T>((uint32_t)m, (uint32_t)g, pass, key, n, 3);
				const int p = mr.part;
				const T xo0 = X[(size_t)p * B + tid], xo1 = X[(size_t)(n + p) * B + tid],
				        xo2 = X[(size_t)(2 * n + p) * B + tid];
				const T xn0 = xo0 + step * mr.z0, xn1 = xo1 + step * mr.z1, xn2 = xo2 + step * mr.z2;
				T d = aP * ((xn0 * xn0 + xn1 * xn1 + xn2 * xn2) - (xo0 * xo0 + xo1 * xo1 + xo2 * xo2));
				for (int i = 0; i < n; i++) {
					const T a0 = X[(size_t)i * B + tid], a1 = X[(size_t)(n + i) * B + tid],
					        a2 = X[(size_t)(2 * n + i) * B + tid];
					const T e0 = a0 - xn0, e1 = a1 - xn1, e2 = a2 - xn2;
					const T f0 = a0 - xo0, f1 = a1 - xo1, f2 = a2 - xo2;
					const T r2n = fma(e2, e2, fma(e1, e1, e0 * e0));
					const T r2o = fma(f2, f2, fma(f1, f1, f0 * f0));
					const T du = drop_u<T>(sy, r2n, coef) - drop_u<T>(sy, r2o, coef);
					d += (i != p) ? du : T(0);
				}
				// exp(2 delta) >= U; a non-finite or overflowing quotient rejects (TDVMC.cpp:886-915)
				const T two = T(2) * d;
				if (isfinite(two) && two >= log(mr.u) && two < (T)kLogDblMax) {
					X[(size_t)p * B + tid] = xn0;
					X[(size_t)(n + p) * B + tid] = xn1;
					X[(size_t)(2 * n + p) * B + tid] = xn2;
					nacc++;
				}
			}
			for (int e = 0; e < 3 * n; e++) pw[e] = X[(size_t)e * B + tid];
			acc_out[g] = nacc;
		}
	}
	(void)nmax;
}

// Cutoff r <= r_max of an FP32 pair decided as FP64 decides it for the same
// coordinates (see within_rmax of the bulk kernels); open boundaries.
template <typename T>
__device__ __forceinline__ bool drop_within(const DropSys& sy, T r, T a0, T a1, T a2, T b0, T b1, T b2) {
	if constexpr (sizeof(T) == 4) {
		if (r > sy.rcut_lo && r < sy.rcut_hi) {
			const double d0 = (double)a0 - (double)b0, d1 = (double)a1 - (double)b1, d2 = (double)a2 - (double)b2;
			return sqrt(fma(d2, d2, fma(d1, d1, d0 * d0))) <= sy.rmax;
		}
	}
	return r <= (T)sy.rmax;
}

// interval and local coordinate on [0, r_max] (uniform knots)
template <typename T>
__device__ __forceinline__ int drop_locate(const DropSys& sy, T r, T& t) {
	if constexpr (sizeof(T) == 4) {
		float jf;
		const int j = floor_clamp(r * sy.hf, sy.nbin - 1, jf);
		t = fmaf(r, sy.hf_lo, fmaf(r, sy.hf, -jf));
		return j;
	} else {
		const T x = r * (T)sy.hinv;
		T jf;
		const int j = floor_clamp(x, sy.nbin - 1, jf);
		t = x - jf;
		return j;
	}
}

// Per-thread shared-memory rows of the evaluation kernel (nmax particles, ns splines,
// ns - 3 knot intervals)
__host__ __device__ inline int drop_eval_rows(int nmax, int ns, bool adj) {
	return 9 * nmax + ns * (adj ? 4 : 1) + 4 * (ns - 3);
}

// Local quantities of every walker of every drop: ln psi, O_k (the folded
// spline sums and O_p = sum |r_i|^2), E_loc, the kinetic sums and, with ADJ,
// dE_loc/d alpha (the same quantities as k_eloc / k_eloc_rev plus the
// one-body and trap terms).  Shared memory: the item's table coefC[nbin_max]
// (three 4-vectors per interval) | rows [drop_eval_rows][blockDim]:
//   X[3 nmax] | G[6 nmax] (gRx gRy gRz gIx gIy gIz per particle) | S[ns] |
//   (ADJ) Lsp[ns] | AR[ns] | AI[ns] | M[4 (ns - 3)]
// M: the forward sweep's moments sum t^c (c = 0..3) of the pairs in each interval,
// turned into the spline sums S and the B'' part of Lsp after the sweep (one
// record update per pair instead of one per spline and sum).
// loc: the uniform piece polynomials [q][c] (also constant for all drops).
template <typename T, bool ADJ>
__global__ void __launch_bounds__(128) k_drop_eval(DropConst dc, const DropSys* __restrict__ sys,
                                                  const int4* __restrict__ items, int nitems,
                                                  int* __restrict__ counter, const T* __restrict__ coefC,
                                                  const double* __restrict__ stage, const double* __restrict__ fold,
                                                  const double* __restrict__ loc, const T* __restrict__ pos, int nmax,
                                                  T* __restrict__ lnpsi_o, T* __restrict__ O_o, T* __restrict__ eloc_o,
                                                  T* __restrict__ other_o, T* __restrict__ dE_o) {
	extern __shared__ __align__(32) unsigned char smem_raw[];
	Q4<T>* cC = reinterpret_cast<Q4<T>*>(smem_raw);
	T* rows = reinterpret_cast<T*>(cC + 3 * dc.nbin_max);
	const int tid = threadIdx.x, B = blockDim.x;
	const int ns = dc.ns, P = dc.p, p1 = dc.p1;
	auto R = [&](int row) -> T& { return rows[(size_t)row * B + tid]; };
	const int oG = 3 * nmax, oS = 9 * nmax, oL = oS + ns, oA = oL + ns, oB = oA + ns;
	const int oM = oS + (ADJ ? 4 : 1) * ns, nbm = ns - 3;
	// uniform pieces: value, first and second derivative in t
	T lv[4][4];
#pragma unroll
	for (int q = 0; q < 4; q++)
#pragma unroll
		for (int c = 0; c < 4; c++) lv[q][c] = (T)loc[q * 4 + c];
	const T dm1 = T(2);
	// the fold's nonzero entries, row by row (a few per row: the boundary rows and
	// one per interior parameter), so each walker's O_k and dE_k sums skip the zeros
	// of the dense [P][ns] matrix; the order of every sum is that of the dense loop
	constexpr int kNnzMax = 4 * (kDropMaxP + 2);
	__shared__ int fk_start[kDropMaxP + 1], fk_sp[kNnzMax];
	__shared__ double fk_f[kNnzMax];
	__shared__ float fk_f32[kNnzMax];
	__shared__ int fk_dense;
	if (tid == 0) {
		int e = 0;
		fk_dense = 0;
		for (int k = 0; k < P; k++) {
			fk_start[k] = e;
			for (int sp = 0; sp < ns; sp++) {
				const double f = fold[(size_t)k * ns + sp];
				if (f == 0.0) continue;
				if (e < kNnzMax) {
					fk_sp[e] = sp;
					fk_f[e] = f;
					fk_f32[e] = (float)f;
				}
				e++;
			}
		}
		fk_start[P] = e;
		fk_dense = e > kNnzMax;
	}
	__syncthreads();
	auto fold_row = [&](int k, int oRow, double scale, int oAdd) -> T {
		// sum over sp of fold[k][sp] * (scale * R(oRow + sp) + R(oAdd + sp)) (oAdd < 0: none),
		// in T: FP32 in the mixed path, the outputs' precision (the FP64 pipe issues a small
		// fraction of the FP32 rate, and the FP64 terms per walker showed in the kernel)
		if constexpr (sizeof(T) == 4) {
			if (!fk_dense) {
				float v = 0.f;
				const float sc = (float)scale;
				for (int e = fk_start[k]; e < fk_start[k + 1]; e++) {
					const int sp = fk_sp[e];
					v += fk_f32[e] * (sc * R(oRow + sp) + (oAdd >= 0 ? R(oAdd + sp) : 0.f));
				}
				return v;
			}
		}
		double v = 0.0;
		if (!fk_dense) {
			for (int e = fk_start[k]; e < fk_start[k + 1]; e++) {
				const int sp = fk_sp[e];
				v += fk_f[e] * (scale * (double)R(oRow + sp) + (oAdd >= 0 ? (double)R(oAdd + sp) : 0.0));
			}
		} else {
			for (int sp = 0; sp < ns; sp++) {
				const double f = fold[(size_t)k * ns + sp];
				if (f == 0.0) continue;
				v += f * (scale * (double)R(oRow + sp) + (oAdd >= 0 ? (double)R(oAdd + sp) : 0.0));
			}
		}
		return (T)v;
	};
	for (;;) {
		const int it = next_item(counter);
		if (it >= nitems) break;
		const int4 wi = items[it];
		const int s = wi.x;
		const DropSys sy = sys[s];
		const int n = sy.n;
		for (int i = tid; i < 3 * sy.nbin; i += B) {
			const T* c = coefC + (size_t)s * dc.nbin_max * 12 + (size_t)i * 4;
			cC[i] = Q4<T>{c[0], c[1], c[2], c[3]};
		}
		const double* prm = stage + (size_t)s * dc.np;
		__syncthreads();
		if (tid >= wi.z) continue;
		const int64_t w = wi.y + tid;
		const int64_t g = (int64_t)s * dc.nws + w;
		const T* pw = pos + sy.pos_off + (size_t)w * 3 * n;
		for (int e = 0; e < 3 * n; e++) R(e) = pw[e];
		for (int e = 0; e < 6 * n; e++) R(oG + e) = T(0);
		for (int k = 0; k < (ADJ ? 4 : 1) * ns; k++) R(oS + k) = T(0);
		for (int k = 0; k < 4 * nbm; k++) R(oM + k) = T(0);
		const T rmaxT = (T)sy.rmax;
		const T hj = (T)sy.hinv;
		KSum<T> vsum, lapR, lapI;
		int nout = 0;
		// forward sweep over unordered pairs (a, i < a); row a's gradient in registers
		for (int a = 1; a < n; a++) {
			const T xa = R(a), ya = R(n + a), za = R(2 * n + a);
			T ga[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
			T lr = T(0), li = T(0), vb = T(0);
			for (int i = 0; i < a; i++) {
				const T xi = R(i), yi = R(n + i), zi = R(2 * n + i);
				const T dx = xa - xi, dy = ya - yi, dz = za - zi;
				const T r2 = fma(dz, dz, fma(dy, dy, dx * dx));
				const T rinv = rsqrt_(r2);
				const T r = r2 * rinv;
				vb += (T)dc.v0 * exp(-r2 * (T)dc.inv2s2);
				if (!drop_within<T>(sy, r, xa, ya, za, xi, yi, zi)) {
					nout++;
					continue;
				}
				T t;
				const int j = drop_locate<T>(sy, r, t);
				const Q4<T> cR = cC[3 * j], cI = cC[3 * j + 1], c2 = cC[3 * j + 2];
				const T d1R = fma(t, fma(t, cR.z, cR.y), cR.x), d1I = fma(t, fma(t, cI.z, cI.y), cI.x);
				const T d2R = fma(t, c2.x, cR.w), d2I = fma(t, c2.y, cI.w);
				const T gR = d1R * rinv, gI = d1I * rinv;
				const T q[6] = {gR * dx, gR * dy, gR * dz, gI * dx, gI * dy, gI * dz};
#pragma unroll
				for (int c = 0; c < 6; c++) {
					ga[c] += q[c];
					R(oG + c * n + i) -= q[c];
				}
				lr += d2R + dm1 * gR;
				li += d2I + dm1 * gI;
				const T t2 = t * t;
				R(oM + 4 * j) += T(1);
				R(oM + 4 * j + 1) += t;
				R(oM + 4 * j + 2) += t2;
				R(oM + 4 * j + 3) += t2 * t;
			}
#pragma unroll
			for (int c = 0; c < 6; c++) R(oG + c * n + a) += ga[c];
			lapR.add(T(2) * lr);
			lapI.add(T(2) * li);
			vsum.add(vb);
		}
		// moments -> spline sums S_s and (ADJ) the B'' part of Lsp: spline s = j + 3 - q on
		// interval j; B'' of both orderings (the (D-1)/r B' part of the Laplacian of O_k enters
		// through the reverse sweep's (D-1)/r term)
		for (int sp = 0; sp < ns; sp++) {
			T sv = T(0), lv2 = T(0);
#pragma unroll
			for (int qq = 0; qq < 4; qq++) {
				const int j = sp - 3 + qq;
				if (j < 0 || j >= nbm) continue;
				const T m0 = R(oM + 4 * j), m1 = R(oM + 4 * j + 1), m2 = R(oM + 4 * j + 2), m3 = R(oM + 4 * j + 3);
				sv += lv[qq][0] * m0 + lv[qq][1] * m1 + lv[qq][2] * m2 + lv[qq][3] * m3;
				if (ADJ) lv2 += T(2) * lv[qq][2] * m0 + T(6) * lv[qq][3] * m1;
			}
			R(oS + sp) = sv;
			if (ADJ) R(oL + sp) = T(2) * hj * hj * lv2;
		}
		// one-body term and trap: gradient 2 alpha_p r, Laplacian 2 D alpha_p per particle
		const T aR = (T)prm[P], aI = (T)prm[p1 + P];
		KSum<T> r2s, e1, e2, e12, gxr, gxi;
		for (int a = 0; a < n; a++) {
			const T x[3] = {R(a), R(n + a), R(2 * n + a)};
			T gr[3], gi[3];
#pragma unroll
			for (int c = 0; c < 3; c++) {
				gr[c] = R(oG + c * n + a) + T(2) * aR * x[c];
				gi[c] = R(oG + (3 + c) * n + a) + T(2) * aI * x[c];
				if (ADJ) {
					R(oG + c * n + a) = gr[c];
					R(oG + (3 + c) * n + a) = gi[c];
				}
			}
			r2s.add(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
			e1.add(gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2]);
			e2.add(gi[0] * gi[0] + gi[1] * gi[1] + gi[2] * gi[2]);
			e12.add(T(2) * (gr[0] * gi[0] + gr[1] * gi[1] + gr[2] * gi[2]));
			gxr.add(gr[0] * x[0] + gr[1] * x[1] + gr[2] * x[2]);
			gxi.add(gi[0] * x[0] + gi[1] * x[1] + gi[2] * x[2]);
		}
		const double c = dc.hbar2_2m;
		const double r2sum = (double)r2s.value();
		const double sR2 = (double)lapR.value() + 6.0 * (double)aR * n;
		const double sI2 = (double)lapI.value() + 6.0 * (double)aI * n;
		const double sR1 = (double)e1.value(), sI1 = (double)e2.value(), sR1I1 = (double)e12.value();
		const double kinR = -(sR1 - sI1 + sR2) * c;
		const double kinI = -(sR1I1 + sI2) * c;
		const double vtot = (double)vsum.value() + dc.kappa * r2sum;
		// O_k: fold of the spline sums (in T, see fold_row), O_p; ln psi in FP64
		double lnp = prm[P - 1] * (double)nout + prm[P] * r2sum;
		for (int k = 0; k < P; k++) {
			const T ok = fold_row(k, oS, 1.0, -1);
			O_o[(size_t)g * p1 + k] = ok;
			lnp += prm[k] * (double)ok;
		}
		O_o[(size_t)g * p1 + P] = (T)r2sum;
		lnpsi_o[g] = (T)lnp;
		eloc_o[2 * g] = (T)(kinR + vtot);
		eloc_o[2 * g + 1] = (T)kinI;
		T* ot = other_o + (size_t)g * 7;
		ot[0] = (T)kinR;
		ot[1] = (T)vtot;
		ot[2] = (T)sR1;
		ot[3] = (T)sI1;
		ot[4] = (T)sR2;
		ot[5] = (T)sI2;
		ot[6] = (T)sR1I1;
		if constexpr (ADJ) {
			// reverse sweep over unordered pairs: sum B'_s(r) ((G_a - G_i) . rhat + (D-1)/r)
			for (int a = 1; a < n; a++) {
				const T xa = R(a), ya = R(n + a), za = R(2 * n + a);
				T ga[6];
#pragma unroll
				for (int cc = 0; cc < 6; cc++) ga[cc] = R(oG + cc * n + a);
				for (int i = 0; i < a; i++) {
					const T xi = R(i), yi = R(n + i), zi = R(2 * n + i);
					const T dx = xa - xi, dy = ya - yi, dz = za - zi;
					const T r2 = fma(dz, dz, fma(dy, dy, dx * dx));
					const T rinv = rsqrt_(r2);
					const T r = r2 * rinv;
					if (!drop_within<T>(sy, r, xa, ya, za, xi, yi, zi)) continue;
					T t;
					const int j = drop_locate<T>(sy, r, t);
					const T gR = ((ga[0] - R(oG + i)) * dx + (ga[1] - R(oG + n + i)) * dy +
					              (ga[2] - R(oG + 2 * n + i)) * dz + dm1) * rinv;
					const T gI = ((ga[3] - R(oG + 3 * n + i)) * dx + (ga[4] - R(oG + 4 * n + i)) * dy +
					              (ga[5] - R(oG + 5 * n + i)) * dz) * rinv;
#pragma unroll
					for (int qq = 0; qq < 4; qq++) {
						const int sp = j + 3 - qq;
						const T b1 = hj * (lv[qq][1] + T(2) * lv[qq][2] * t + T(3) * lv[qq][3] * t * t);
						R(oA + sp) += b1 * gR;
						R(oB + sp) += b1 * gI;
					}
				}
			}
			for (int k = 0; k < P; k++) {
				const T re = fold_row(k, oA, 2.0, oL), im = fold_row(k, oB, 2.0, -1);
				dE_o[((size_t)g * p1 + k) * 2 + 0] = (T)(-c) * re;
				dE_o[((size_t)g * p1 + k) * 2 + 1] = (T)(-c) * im;
			}
			dE_o[((size_t)g * p1 + P) * 2 + 0] = (T)(-c * (6.0 * n + 4.0 * (double)gxr.value()));
			dE_o[((size_t)g * p1 + P) * 2 + 1] = (T)(-c * 4.0 * (double)gxi.value());
		}
	}
}

// Per-drop walker means and centred second moments (one block per drop):
// pass 1 the means of the DropCols columns (FP64 sums in a fixed order; FP32
// inputs summed per chunk with carried rounding errors), pass 2
// S_kl = <(O_k - <O_k>)(O_l - <O_l>)> and cov(O_k, E^R), cov(O_k, E^I).  The
// centred products are formed in T and summed in T over runs of 32 walkers,
// each run added in FP64 (FP64 issue is scarce on this GPU).  Both passes stage
// the drop's walkers in chunks of kDropRedStage through shared memory: each
// per-walker array (O, E, the other values, the acceptance count, dE) is one
// contiguous range of global memory for a chunk, copied as such (coalesced,
// several loads in flight per thread, no per-element column arithmetic), and a
// summing thread reads its column with a fixed base and stride.  The order of
// every sum is that of a walker-by-walker loop.
constexpr int kDropReduceThreads = 256;
constexpr int kDropRedChunk = 32;   // walkers per pass-2 run
constexpr int kDropRedStage = 128;  // walkers per staged chunk (whole runs)
constexpr int kDropCols = 3 * (kDropMaxP + 1) + 10;   // DropCols count at the largest p
constexpr int kDropEntries = (kDropMaxP + 1) * (kDropMaxP + 2) / 2 + 2 * (kDropMaxP + 1);
constexpr int kDropEntriesPerThread = (kDropEntries + kDropReduceThreads - 1) / kDropReduceThreads;
// pass 1: the four interleaved partial sums of a column (walkers w = q mod 4) are
// summed by four threads
constexpr int kDropMeanSlots = (4 * kDropCols + kDropReduceThreads - 1) / kDropReduceThreads;
static_assert(kDropRedStage % 4 == 0 && kDropRedStage % kDropRedChunk == 0, "chunks of whole runs and phases");

// dst[0, count) <- src[0, count) by the block's threads
template <typename D, typename S>
__device__ __forceinline__ void red_copy(D* __restrict__ dst, const S* __restrict__ src, int count, int tid) {
#pragma unroll 4
	for (int e = tid; e < count; e += kDropReduceThreads) dst[e] = (D)src[e];
}

template <typename T>
__global__ void __launch_bounds__(kDropReduceThreads) k_drop_reduce(
    DropConst dc, const T* __restrict__ O, const T* __restrict__ eloc, const T* __restrict__ other7,
    const int* __restrict__ acc, const T* __restrict__ dE, int use_dE, double* __restrict__ means,
    double* __restrict__ S, double* __restrict__ cov) {
	__shared__ double m_s[kDropCols];
	__shared__ double part_s[4 * kDropCols];
	// staged chunk: sO[cw p1] | sE[2 cw] | sX[7 cw] | sA[cw] | sD[2 p1 cw]
	extern __shared__ __align__(16) unsigned char red_raw[];
	const int s = blockIdx.x, tid = threadIdx.x;
	const int p1 = dc.p1;
	const DropCols cl{p1};
	const int K = cl.count();
	T* sO = reinterpret_cast<T*>(red_raw);
	T* sE = sO + (size_t)kDropRedStage * p1;
	T* sX = sE + 2 * kDropRedStage;
	T* sA = sX + 7 * kDropRedStage;
	T* sD = sA + kDropRedStage;
	const int64_t g0 = (int64_t)s * dc.nws, nw = dc.nws;
	// pass 1: slot (column c, phase q) sums walkers w = q mod 4 of column c in FP64,
	// the four interleaved sums of a walker-by-walker loop; a thread owns
	// kDropMeanSlots slots (tid + k blockDim)
	const T* cb[kDropMeanSlots];  // the slot's column: cb[w * cs]
	int cs[kDropMeanSlots], cq[kDropMeanSlots];
	bool live[kDropMeanSlots];
	double a[kDropMeanSlots];
#pragma unroll
	for (int k = 0; k < kDropMeanSlots; k++) {
		const int slot = tid + k * kDropReduceThreads, c = slot >> 2;
		cq[k] = slot & 3;
		a[k] = 0.0;
		cb[k] = sO;
		cs[k] = 0;
		live[k] = c < K;
		if (c < p1) {
			cb[k] = sO + c;
			cs[k] = p1;
		} else if (c < cl.other()) {
			cb[k] = sE + (c - cl.ER());
			cs[k] = 2;
		} else if (c < cl.acc()) {
			cb[k] = sX + (c - cl.other());
			cs[k] = 7;
		} else if (c == cl.acc()) {
			cb[k] = sA;
			cs[k] = 1;
		} else if (c < K) {
			cb[k] = sD + (c - cl.dE());
			cs[k] = 2 * p1;
			live[k] = use_dE != 0;
		}
	}
	for (int64_t w0 = 0; w0 < nw; w0 += kDropRedStage) {
		const int cw = (int)(nw - w0 < kDropRedStage ? nw - w0 : kDropRedStage);
		const int64_t g = g0 + w0;
		__syncthreads();
		red_copy(sO, O + (size_t)g * p1, cw * p1, tid);
		red_copy(sE, eloc + 2 * (size_t)g, 2 * cw, tid);
		red_copy(sX, other7 + 7 * (size_t)g, 7 * cw, tid);
		red_copy(sA, acc + g, cw, tid);
		if (use_dE) red_copy(sD, dE + (size_t)g * 2 * p1, 2 * p1 * cw, tid);
		__syncthreads();
		// w0 is a multiple of 4, so walker w of the chunk has phase w mod 4.  FP32: the
		// slot's walkers of the chunk are summed in FP32 with the error of every addition
		// carried (two-sum), and the chunk's sum and error are added in FP64 (with one FP64
		// addition per walker, FP64 issue bounded the pass: 0.71 -> 0.37 ms per stage)
#pragma unroll
		for (int k = 0; k < kDropMeanSlots; k++) {
			if (!live[k]) continue;
			if constexpr (sizeof(T) == 4) {
				float sum = 0.f, err = 0.f;
				for (int w = cq[k]; w < cw; w += 4) {
					const float x = cb[k][(size_t)w * cs[k]];
					const float t = sum + x, bp = t - sum;
					err += (sum - (t - bp)) + (x - bp);
					sum = t;
				}
				a[k] += (double)sum + (double)err;
			} else {
				for (int w = cq[k]; w < cw; w += 4) a[k] += (double)cb[k][(size_t)w * cs[k]];
			}
		}
	}
#pragma unroll
	for (int k = 0; k < kDropMeanSlots; k++) {
		const int slot = tid + k * kDropReduceThreads;
		if (slot < 4 * K) part_s[slot] = a[k];
	}
	__syncthreads();
	if (tid < K) {
		const double* pq = part_s + 4 * tid;
		const double mval = ((pq[0] + pq[1]) + (pq[2] + pq[3])) / (double)nw;
		m_s[tid] = mval;
		means[(size_t)s * K + tid] = mval;
	}
	__syncthreads();
	// pass 2: thread per entry of the upper triangle of S and the two covariance
	// columns (column p1: E^R, p1 + 1: E^I), each factor centred in T as it is read
	const int nS = p1 * (p1 + 1) / 2, nE = nS + 2 * p1;
	const T* bi[kDropEntriesPerThread];
	const T* bj[kDropEntriesPerThread];
	int si[kDropEntriesPerThread], sj[kDropEntriesPerThread], ei[kDropEntriesPerThread], ej[kDropEntriesPerThread];
	T mi[kDropEntriesPerThread], mj[kDropEntriesPerThread];
	double acc64[kDropEntriesPerThread];
#pragma unroll
	for (int q = 0; q < kDropEntriesPerThread; q++) {
		const int e = tid + q * kDropReduceThreads;
		int i = 0, j = 0;
		if (e < nS) {
			// row-major upper triangle: e -> (i, j), j >= i
			int rem = e;
			while (rem >= p1 - i) {
				rem -= p1 - i;
				i++;
			}
			j = i + rem;
		} else if (e < nE) {
			i = (e - nS) >> 1;
			j = p1 + ((e - nS) & 1);
		}
		ei[q] = i;
		ej[q] = j;
		bi[q] = sO + i;
		si[q] = p1;
		mi[q] = (T)m_s[i];
		if (j < p1) {
			bj[q] = sO + j;
			sj[q] = p1;
			mj[q] = (T)m_s[j];
		} else {
			bj[q] = sE + (j - p1);
			sj[q] = 2;
			mj[q] = (T)m_s[j == p1 ? cl.ER() : cl.EI()];
		}
		acc64[q] = 0.0;
	}
	for (int64_t w0 = 0; w0 < nw; w0 += kDropRedStage) {
		const int cw = (int)(nw - w0 < kDropRedStage ? nw - w0 : kDropRedStage);
		const int64_t g = g0 + w0;
		__syncthreads();
		red_copy(sO, O + (size_t)g * p1, cw * p1, tid);
		red_copy(sE, eloc + 2 * (size_t)g, 2 * cw, tid);
		__syncthreads();
		// runs of kDropRedChunk walkers in order, each summed in T and added in FP64
		for (int r0 = 0; r0 < cw; r0 += kDropRedChunk) {
			const int r1 = r0 + kDropRedChunk < cw ? r0 + kDropRedChunk : cw;
#pragma unroll
			for (int q = 0; q < kDropEntriesPerThread; q++) {
				if (tid + q * kDropReduceThreads >= nE) break;
				T run = T(0);
				for (int w = r0; w < r1; w++)
					run = fma(bi[q][(size_t)w * si[q]] - mi[q], bj[q][(size_t)w * sj[q]] - mj[q], run);
				acc64[q] += (double)run;
			}
		}
	}
#pragma unroll
	for (int q = 0; q < kDropEntriesPerThread; q++) {
		const int e = tid + q * kDropReduceThreads;
		if (e >= nE) break;
		const double v = acc64[q] / (double)nw;
		if (e < nS) {
			S[(size_t)s * p1 * p1 + (size_t)ei[q] * p1 + ej[q]] = v;
			S[(size_t)s * p1 * p1 + (size_t)ej[q] * p1 + ei[q]] = v;
		} else {
			cov[((size_t)s * p1 + ei[q]) * 2 + (ej[q] - p1)] = v;
		}
	}
}

}  // namespace tdvmc
