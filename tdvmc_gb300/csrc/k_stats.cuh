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

// Column col of walker w in the pass-1 layout (the wf column, exp(ln psi + phi^R),
// comes from wfv: the block's exponentials, computed lane-parallel beforehand
// because FP64 issue is scarce and exp is dozens of FP64 instructions).
template <typename T>
__device__ __forceinline__ T cols1_value(const Cols1& c, int col, int64_t w, const T* __restrict__ O,
                                         const T* __restrict__ eloc, const T* __restrict__ other7,
                                         const T* __restrict__ lnpsi, const int* __restrict__ acc,
                                         const T* __restrict__ dE, int use_dE) {
	const int p = c.p;
	if (col < p) return O[(size_t)w * p + col];
	if (col == c.ER()) return eloc[2 * w];
	if (col == c.EI()) return eloc[2 * w + 1];
	if (col < c.wf()) return other7[(size_t)w * 7 + (col - c.other())];
	if (col == c.lnpsi()) return lnpsi[w];
	if (col == c.acc()) return (T)acc[w];
	return use_dE ? dE[(size_t)w * 2 * p + (col - c.dE())] : T(0);
}

// Pass 1: one thread per column over the block's walker range, four
// independent FP64 running sums added in a fixed order (every walker's value
// enters an FP64 sum directly, so FP32 inputs are added without FP32 rounding).
constexpr int kReduce1MaxWalkers = 64;  // walkers per block (shared exponentials)
template <typename T>
__global__ void __launch_bounds__(256) k_reduce1(int p, int64_t nw, const T* __restrict__ O, const T* __restrict__ eloc,
                                                 const T* __restrict__ other7, const T* __restrict__ lnpsi,
                                                 const int* __restrict__ acc, const T* __restrict__ dE, int use_dE,
                                                 const double* __restrict__ params, double* __restrict__ partial) {
	__shared__ double wfv[kReduce1MaxWalkers];
	Cols1 c{p};
	const int K = c.count();
	const int64_t per = (nw + gridDim.x - 1) / gridDim.x;
	const int64_t w0 = (int64_t)blockIdx.x * per;
	const int64_t w1 = (w0 + per < nw) ? w0 + per : nw;
	const double phiR = params[2 * p];
	const int nloc = (int)(w1 > w0 ? w1 - w0 : 0);
	for (int i = threadIdx.x; i < nloc; i += blockDim.x) wfv[i] = exp((double)lnpsi[w0 + i] + phiR);
	__syncthreads();
	for (int col = threadIdx.x; col < K; col += blockDim.x) {
		double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
		if (col == c.wf()) {
			int i = 0;
			for (; i + 4 <= nloc; i += 4) {
				s0 += wfv[i];
				s1 += wfv[i + 1];
				s2 += wfv[i + 2];
				s3 += wfv[i + 3];
			}
			for (; i < nloc; i++) s0 += wfv[i];
		} else {
			int64_t w = w0;
			for (; w + 4 <= w1; w += 4) {
				s0 += (double)cols1_value(c, col, w, O, eloc, other7, lnpsi, acc, dE, use_dE);
				s1 += (double)cols1_value(c, col, w + 1, O, eloc, other7, lnpsi, acc, dE, use_dE);
				s2 += (double)cols1_value(c, col, w + 2, O, eloc, other7, lnpsi, acc, dE, use_dE);
				s3 += (double)cols1_value(c, col, w + 3, O, eloc, other7, lnpsi, acc, dE, use_dE);
			}
			for (; w < w1; w++) s0 += (double)cols1_value(c, col, w, O, eloc, other7, lnpsi, acc, dE, use_dE);
		}
		partial[(size_t)blockIdx.x * K + col] = (s0 + s1) + (s2 + s3);
	}
}

// Sum `nblk` partial rows of width K in fixed order and scale by `scale`: one
// warp per column, lane l adding rows l, l + 32, ..., then a fixed butterfly.
constexpr int kFinalizeThreads = 256;
__global__ void __launch_bounds__(kFinalizeThreads) k_finalize(int K, int nblk, const double* __restrict__ partial,
                                                               double scale, double* __restrict__ out) {
	const int lane = threadIdx.x & 31;
	const int col = blockIdx.x * (kFinalizeThreads / 32) + (threadIdx.x >> 5);
	if (col >= K) return;  // whole warps
	double s = 0.0;
	for (int b = lane; b < nblk; b += 32) s += partial[(size_t)b * K + col];
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
	if (lane == 0) out[col] = s * scale;
}
inline int finalize_blocks(int K) { return (K + kFinalizeThreads / 32 - 1) / (kFinalizeThreads / 32); }

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
	if (with_S) {
		for (int e = threadIdx.x; e < npair; e += blockDim.x) {
			const int k = e / ncol, l = e % ncol;
			double s = 0.0;
			for (int r = 0; r < nt; r++) s += ytile[r * ncol + k] * ytile[r * ncol + l];
			partial[(size_t)blockIdx.x * npair + e] = s;
		}
		return;
	}
	// only the energy columns l = p, p + 1; four lanes per entry (rows r = q mod 4),
	// added in a fixed order; the S block of the row stays zero
	for (int e = threadIdx.x; e < npair; e += blockDim.x)
		if (e % ncol < p) partial[(size_t)blockIdx.x * npair + e] = 0.0;
	for (int t = threadIdx.x; t < ((2 * p * 4 + 31) & ~31); t += blockDim.x) {
		const int e2 = t >> 2, q = t & 3;
		const bool on = e2 < 2 * p;
		const int k = on ? e2 >> 1 : 0, l = p + (e2 & 1);
		double s = 0.0;
		if (on)
			for (int r = q; r < nt; r += 4) s += ytile[r * ncol + k] * ytile[r * ncol + l];
		s += __shfl_xor_sync(0xffffffffu, s, 1);
		s += __shfl_xor_sync(0xffffffffu, s, 2);
		if (on && q == 0) partial[(size_t)blockIdx.x * npair + k * ncol + l] = s;
	}
}

}  // namespace tdvmc
