// Walker-mean statistics: the single-GPU replacement of the per-rank
// accumulation (UpdateExpectationValues, TDVMC.cpp:1103-1109) plus the MPI
// ReduceToAverage (TDVMC.cpp:1182-1188, MPIMethods.h:191-206).
//
// Two deterministic passes, each a grid of blocks writing FP64 partial sums
// followed by one block that adds the partials in fixed order:
//   pass 1  means of O_k, E^R, E^I, the kinetic partial sums, wf, ln psi,
//           the acceptance count and (adjoint) dE_loc/d alpha;
//   pass 2  centred second moments: S_kl = <(O_k - <O_k>)(O_l - <O_l>)> and
//           the covariances of O_k with E^R and E^I, in FP64.
// The mixed-precision path replaces the S block of pass 2 by the 3xTF32
// tensor-core contraction of k_gram_tf32.cuh; the covariances stay FP64.
#pragma once

#include "common.cuh"

namespace tdvmc {

// Column layout of pass 1 (K1 = 3p + 12 columns).
struct Cols1 {
	int p;
	__host__ __device__ int O() const { return 0; }
	__host__ __device__ int ER() const { return p; }
	__host__ __device__ int EI() const { return p + 1; }
	__host__ __device__ int other() const { return p + 2; }  // 7
	__host__ __device__ int wf() const { return p + 9; }
	__host__ __device__ int lnpsi() const { return p + 10; }
	__host__ __device__ int acc() const { return p + 11; }
	__host__ __device__ int dE() const { return p + 12; }  // 2p
	__host__ __device__ int count() const { return 3 * p + 12; }
};

template <typename T>
__global__ void __launch_bounds__(256) k_reduce1(int p, int64_t nw, const T* __restrict__ O, const T* __restrict__ eloc,
                                                 const T* __restrict__ other7, const T* __restrict__ lnpsi,
                                                 const int* __restrict__ acc, const T* __restrict__ dE, int use_dE,
                                                 const double* __restrict__ params, double* __restrict__ partial) {
	Cols1 c{p};
	const int K = c.count();
	const int64_t per = (nw + gridDim.x - 1) / gridDim.x;
	const int64_t w0 = (int64_t)blockIdx.x * per;
	const int64_t w1 = (w0 + per < nw) ? w0 + per : nw;
	const double phiR = params[2 * p];
	for (int col = threadIdx.x; col < K; col += blockDim.x) {
		double s = 0.0;
		for (int64_t w = w0; w < w1; w++) {
			double v;
			if (col < p) v = (double)O[(size_t)w * p + col];
			else if (col == c.ER()) v = (double)eloc[2 * w];
			else if (col == c.EI()) v = (double)eloc[2 * w + 1];
			else if (col < c.wf()) v = (double)other7[(size_t)w * 7 + (col - c.other())];
			else if (col == c.wf()) v = exp((double)lnpsi[w] + phiR);
			else if (col == c.lnpsi()) v = (double)lnpsi[w];
			else if (col == c.acc()) v = (double)acc[w];
			else v = use_dE ? (double)dE[(size_t)w * 2 * p + (col - c.dE())] : 0.0;
			s += v;
		}
		partial[(size_t)blockIdx.x * K + col] = s;
	}
}

// Sum `nblk` partial rows of width K in fixed order and scale by `scale`.
__global__ void __launch_bounds__(256) k_finalize(int K, int nblk, const double* __restrict__ partial, double scale,
                                                  double* __restrict__ out) {
	for (int col = threadIdx.x; col < K; col += blockDim.x) {
		double s = 0.0;
		for (int b = 0; b < nblk; b++) s += partial[(size_t)b * K + col];
		out[col] = s * scale;
	}
}

// Pass 2 (FP64): Y = [O - <O> | E^R - <E^R> | E^I - <E^I>] (p + 2 columns).
// Block b stages walkers [b*chunk, (b+1)*chunk) of Y in shared memory and
// writes partial[b] = (Y^T Y)[0..p-1][0..p+1] (with_S = 0: only the two
// energy columns, the S block being computed elsewhere).
template <typename T>
__global__ void __launch_bounds__(256) k_reduce2(int p, int64_t nw, int chunk, const T* __restrict__ O,
                                                 const T* __restrict__ eloc, const double* __restrict__ means,
                                                 int with_S, double* __restrict__ partial) {
	extern __shared__ double ytile[];  // [chunk][p + 2]
	const int ncol = p + 2;
	const int64_t w0 = (int64_t)blockIdx.x * chunk;
	const int nt = (int)((nw - w0) < chunk ? (nw - w0) : chunk);
	for (int e = threadIdx.x; e < nt * ncol; e += blockDim.x) {
		const int r = e / ncol, col = e % ncol;
		const int64_t w = w0 + r;
		double v;
		if (col < p) v = (double)O[(size_t)w * p + col] - means[col];
		else if (col == p) v = (double)eloc[2 * w] - means[p];
		else v = (double)eloc[2 * w + 1] - means[p + 1];
		ytile[r * ncol + col] = v;
	}
	__syncthreads();
	const int npair = p * ncol;
	for (int e = threadIdx.x; e < npair; e += blockDim.x) {
		const int k = e / ncol, l = e % ncol;
		double s = 0.0;
		if (with_S || l >= p)
			for (int r = 0; r < nt; r++) s += ytile[r * ncol + k] * ytile[r * ncol + l];
		partial[(size_t)blockIdx.x * npair + e] = s;
	}
}

}  // namespace tdvmc
