// Walker statistics for callers that cannot allocate device memory.
//
// Some host programs own every byte of GPU memory through their own pool
// allocator and forbid cudaMalloc / cudaFree while they run: a solver
// framework that hands this library slices of its pool, or an embedding
// that must not change the device's memory footprint after start-up.  Such a
// caller can still pass device arrays it already owns.  This entry point
// computes the same FP64 walker means, centred S and energy covariances as
// tdvmc_reduce_stats from caller-owned device arrays, and keeps its per-block
// partial sums in one fixed, file-scope device array instead of allocating.
//
// The array holds kNaScratch doubles (about 0.6 MB) on every device that
// loads this library, until the process exits.  Every call shares it: a
// block writes (not adds) each of its partial sums before they are read, so
// nothing has to start at zero, but two calls whose kernels overlap on the
// GPU (different streams, or different host threads) race on it.
#include "../../include/tdvmc_gpu.h"

#include <cuda_runtime.h>

#include <mutex>

namespace {

constexpr int kNaMaxP = 32;                    // parameters supported
constexpr int kNaCols = kNaMaxP + 2;           // O_k, E^R, E^I
constexpr int kNaBlocks = 64;                  // walker chunks (partial sums)
constexpr int kNaTile = 64;                    // walkers staged per pass-2 tile
constexpr size_t kNaPass1 = (size_t)kNaBlocks * kNaCols;
constexpr size_t kNaScratch = kNaPass1 + (size_t)kNaBlocks * kNaMaxP * kNaCols;

__device__ __align__(256) double g_na_scratch[kNaScratch];

// device address of g_na_scratch per device, looked up once with that device current
constexpr int kNaMaxDevices = 64;
double* g_na_addr[kNaMaxDevices] = {nullptr};
std::mutex g_na_mutex;

__global__ void __launch_bounds__(256) na_pass1(const double* __restrict__ O, const double* __restrict__ eloc,
                                                int64_t nw, int p, int64_t chunk, double* __restrict__ part) {
	const int ncol = p + 2;
	const int64_t w0 = (int64_t)blockIdx.x * chunk;
	const int64_t w1 = (w0 + chunk < nw) ? w0 + chunk : nw;
	for (int c = threadIdx.x; c < ncol; c += blockDim.x) {
		double s = 0.0;
		for (int64_t w = w0; w < w1; w++) s += (c < p) ? O[(size_t)w * p + c] : eloc[2 * w + (c - p)];
		part[(size_t)blockIdx.x * ncol + c] = s;
	}
}

__global__ void __launch_bounds__(256) na_means(int p, int nblk, int64_t nw, const double* __restrict__ part,
                                                double* __restrict__ O_mean, double* __restrict__ E_mean) {
	const int ncol = p + 2;
	for (int c = threadIdx.x; c < ncol; c += blockDim.x) {
		double s = 0.0;
		for (int b = 0; b < nblk; b++) s += part[(size_t)b * ncol + c];
		s /= (double)nw;
		if (c < p) O_mean[c] = s;
		else E_mean[c - p] = s;
	}
}

__global__ void __launch_bounds__(256) na_pass2(const double* __restrict__ O, const double* __restrict__ eloc,
                                                int64_t nw, int p, int64_t chunk, const double* __restrict__ O_mean,
                                                const double* __restrict__ E_mean, double* __restrict__ part) {
	__shared__ double y[kNaTile * kNaCols];
	const int ncol = p + 2;
	const int npair = p * ncol;
	const int64_t w0 = (int64_t)blockIdx.x * chunk;
	const int64_t w1 = (w0 + chunk < nw) ? w0 + chunk : nw;
	double acc[(kNaMaxP * kNaCols + 255) / 256];
#pragma unroll
	for (int q = 0; q < (kNaMaxP * kNaCols + 255) / 256; q++) acc[q] = 0.0;
	for (int64_t tb = w0; tb < w1; tb += kNaTile) {
		const int nt = (int)((w1 - tb) < kNaTile ? (w1 - tb) : kNaTile);
		for (int e = threadIdx.x; e < nt * ncol; e += blockDim.x) {
			const int r = e / ncol, c = e % ncol;
			const int64_t w = tb + r;
			y[r * ncol + c] = (c < p) ? O[(size_t)w * p + c] - O_mean[c] : eloc[2 * w + (c - p)] - E_mean[c - p];
		}
		__syncthreads();
#pragma unroll
		for (int q = 0; q < (kNaMaxP * kNaCols + 255) / 256; q++) {
			const int e = threadIdx.x + q * 256;
			if (e < npair) {
				const int k = e / ncol, l = e % ncol;
				double s = 0.0;
				for (int r = 0; r < nt; r++) s += y[r * ncol + k] * y[r * ncol + l];
				acc[q] += s;
			}
		}
		__syncthreads();
	}
#pragma unroll
	for (int q = 0; q < (kNaMaxP * kNaCols + 255) / 256; q++) {
		const int e = threadIdx.x + q * 256;
		if (e < npair) part[(size_t)blockIdx.x * npair + e] = acc[q];
	}
}

__global__ void __launch_bounds__(256) na_cov(int p, int nblk, int64_t nw, const double* __restrict__ part,
                                              double* __restrict__ S, double* __restrict__ cov_OER,
                                              double* __restrict__ cov_OEI) {
	const int ncol = p + 2;
	const int npair = p * ncol;
	for (int e = threadIdx.x; e < npair; e += blockDim.x) {
		double s = 0.0;
		for (int b = 0; b < nblk; b++) s += part[(size_t)b * npair + e];
		s /= (double)nw;
		const int k = e / ncol, l = e % ncol;
		if (l < p) S[(size_t)k * p + l] = s;
		else if (l == p) cov_OER[k] = s;
		else cov_OEI[k] = s;
	}
}

}  // namespace

extern "C" int tdvmc_reduce_walkers_noalloc(const double* O, const double* eloc, int64_t nw, int32_t p,
                                            double* O_mean, double* E_mean, double* S, double* cov_OER,
                                            double* cov_OEI, void* stream) {
	if (!O || !eloc || !O_mean || !E_mean || !S || !cov_OER || !cov_OEI) return TDVMC_ERR_ARG;
	if (p < 1 || p > kNaMaxP || nw < 1) return TDVMC_ERR_ARG;
	// an error left by the caller's own earlier CUDA work is not this call's:
	// report it without launching and without clearing it
	if (cudaPeekAtLastError() != cudaSuccess) return TDVMC_ERR_CUDA;
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) return TDVMC_ERR_CUDA;
	double* scratch = nullptr;
	{
		std::lock_guard<std::mutex> lock(g_na_mutex);
		if (!g_na_addr[dev]) {
			// a host-side name of a __device__ array is not a device address:
			// look the address up once per device, with that device current
			void* ptr = nullptr;
			if (cudaGetSymbolAddress(&ptr, g_na_scratch) != cudaSuccess || !ptr) return TDVMC_ERR_CUDA;
			g_na_addr[dev] = static_cast<double*>(ptr);
		}
		scratch = g_na_addr[dev];
	}
	cudaStream_t st = static_cast<cudaStream_t>(stream);
	const int nblk = (int)(nw < kNaBlocks ? nw : kNaBlocks);
	const int64_t chunk = (nw + nblk - 1) / nblk;
	double* part1 = scratch;
	double* part2 = scratch + kNaPass1;
	na_pass1<<<nblk, 256, 0, st>>>(O, eloc, nw, p, chunk, part1);
	na_means<<<1, 256, 0, st>>>(p, nblk, nw, part1, O_mean, E_mean);
	na_pass2<<<nblk, 256, 0, st>>>(O, eloc, nw, p, chunk, O_mean, E_mean, part2);
	na_cov<<<1, 256, 0, st>>>(p, nblk, nw, part2, S, cov_OER, cov_OEI);
	return cudaGetLastError() == cudaSuccess ? TDVMC_OK : TDVMC_ERR_CUDA;
}
